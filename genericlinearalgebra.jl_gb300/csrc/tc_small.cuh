// Double-float products of the batched refinement (n <= 128) on the tcgen05
// tensor cores, run by the whole CTA that refines the matrix (no counterpart
// in GenericLinearAlgebra.jl).
//
//   C = P Q,  P (n x n) and Q (n x n) read through accessors returning float
//   pairs, C handed to a store functor as float pairs,
//
// by the Ozaki scheme of the large path's GEMM (ozaki.cuh; K. Ozaki,
// T. Ogita, S. Oishi, S. M. Rump, Numer. Algorithms 59 (2012)): every row i
// of P is scaled by 2^e_i >= max_k |p_ik| and every column j of Q by
// 2^f_j >= max_k |q_kj|, each scaled value is split into seven 7-bit integer
// slices (exact in bf16), and the 28 slice pairs with s + t <= 8 are
// multiplied by tcgen05.mma kind::f16 (bf16 in, FP32 out) into seven "level"
// accumulators in TMEM, L = s + t, each an exact integer sum (K <= 128: at
// most 128 x 37,895 < 2^24, see ozaki.cuh). C_ij = 2^(e_i + f_j) sum_L
// level_L(i, j) 2^(-7 L), summed in double-float: ~2^-47 relative to
// max_k |p_ik| max_k |q_kj| per term, as the double-float SIMT products.
//
// Shape: M = 128 rows of C per MMA (rows >= n are zero slices), N = 32
// columns per pass (7 levels x 32 = 224 of the CTA's 256 TMEM columns; two
// CTAs per SM share the 512), K in slabs of 32. Per pass and slab the CTA
// slices P's 128 x 32 block and Q's 32 x 32 block into shared memory in the
// MMA's canonical no-swizzle K-major layout (oz_prims.cuh), one thread
// issues the MMAs (per K = 16 step one per slice of P, see idesc_n) and
// commits to an mbarrier, and the CTA loads the next slab's values into
// registers while they run; after the last slab the eight warps drain the
// levels with tcgen05.ld (warp w reads TMEM lanes 32 (w % 4) .. +31,
// columns 16 (w / 4) .. +15), combine them and call the store functor.
// With a per-CTA global scratch (the persistent kernel), P's slabs are
// sliced only in the first pass and stored there by bulk copies; later
// passes bring them back with bulk copies and slice only Q's slab.
//
// Every mbarrier wait is bounded: a wait that runs out sets the error word
// and the CTA's abort flag, no further MMA is issued by the CTA, and the
// caller sees `false` (the matrix is then reported as not converged).
// teardown() waits (bounded) for every bulk copy and MMA the CTA issued
// before it frees the TMEM.
#pragma once
#include <cuda_bf16.h>

#include "df64.cuh"
#include "oz_prims.cuh"

namespace gla {
namespace tcs {

constexpr int kS = 7;                       // slices per operand
constexpr int kM = 128;                     // MMA M (rows of C per pass)
constexpr int kNT = 32;                     // columns of C per pass
constexpr int kTmemCols = 256;              // per CTA (two CTAs per SM)
constexpr int kKS = oz::kKS;                // k per slab
constexpr int kABlk = kM * kKS * 2;         // one slice of a P slab: 8 KB
constexpr int kBBlk = kNT * kKS * 2;        // one slice of a Q slab: 2 KB
constexpr int kSmem = kS * (kABlk + kBBlk);  // 70 KB of dynamic shared memory
// kind::f16 instruction descriptor: F32 accumulate (bit 4), bf16 A and B
// (bits 7, 10), both K-major, N >> 3 at bit 17, M >> 4 at bit 24. One MMA
// per A slice s multiplies it by Q's slices 1 .. 8 - s at once: those are
// adjacent 32-row blocks in shared memory (one operand of N = 32 (8 - s)
// rows in the same canonical layout) and their levels s + 1 .. 8 are
// adjacent 32-column accumulators in TMEM.
GLA_DEV constexpr uint32_t idesc_n(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kM >> 4) << 24);
}
static_assert(kS * kNT <= kTmemCols, "level accumulators exceed the CTA's TMEM columns");
// Per-CTA global scratch of P's slices (all slabs of an order-128 operand):
// pass 0 slices P and stores each slab's slices there with a bulk copy;
// later passes load them back with a bulk copy instead of slicing again.
constexpr int kPSlab = kS * kABlk;                 // 56 KB: P's part of a slab
constexpr int kPCacheBytes = (128 / kKS) * kPSlab;  // 224 KB per CTA
static_assert(kM <= 128, "one row of C per TMEM lane");

// Per-CTA state in static shared memory.
struct Shared {
  uint64_t bar;  // MMA completion (one phase per commit)
  uint64_t fin;  // teardown: every MMA of the CTA finished
  uint64_t ldbar;  // bulk loads of cached P slabs (one phase per load)
  uint32_t tmem;
  int abort;
  int ld_pending;  // a bulk load whose completion was not seen (abort path)
  uint32_t ld_parity;
};

struct Ctx {
  Shared* sh;
  unsigned char* slabs;  // kSmem bytes of dynamic shared memory, 16-byte aligned
  unsigned char* pcache; // kPCacheBytes of global scratch of this CTA, or null (no P cache)
  int* err;              // error word in global memory
  uint32_t phase;        // parity of the next completion of sh->bar
  uint32_t ldphase;      // parity of the next completion of sh->ldbar
};

GLA_DEV void bulk_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(oz::smem_u32(ssrc)),
               "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
// the bulk stores of this thread have read their shared-memory source
GLA_DEV void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// the bulk stores of this thread are complete
GLA_DEV void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// All threads of the CTA (256); TMEM is held until teardown().
GLA_DEV void setup(Ctx& c, Shared* sh, unsigned char* slabs, int* err, unsigned char* pcache = nullptr) {
  c.sh = sh;
  c.slabs = slabs;
  c.pcache = pcache;
  c.err = err;
  c.phase = 0;
  c.ldphase = 0;
  if (threadIdx.x == 0) {
    oz::mbar_init(&sh->bar, 1);
    oz::mbar_init(&sh->fin, 1);
    oz::mbar_init(&sh->ldbar, 1);
    sh->abort = 0;
    sh->ld_pending = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(oz::smem_u32(&sh->tmem)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
}

// All threads of the CTA, once, before it exits.
GLA_DEV void teardown(Ctx& c) {
  __syncthreads();
  if (threadIdx.x == 0) {  // the thread that issued every MMA and bulk copy of this CTA
    bulk_wait_all();
    if (c.sh->ld_pending)  // (abort path) the last bulk load lands before the CTA exits
      for (long long it = 0; it < oz::kWaitLimit && !oz::mbar_try(&c.sh->ldbar, c.sh->ld_parity); it++) {
      }
    oz::mma_commit(&c.sh->fin);
    for (long long it = 0; it < oz::kWaitLimit && !oz::mbar_try(&c.sh->fin, 0); it++) {
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(c.sh->tmem), "r"(kTmemCols));
}

GLA_DEV bool ok(const Ctx& c) { return !c.sh->abort; }

// Wait for the next commit (all threads); false once the CTA has aborted.
GLA_DEV bool wait_mma(Ctx& c) {
  if (!c.sh->abort && !oz::mbar_wait(&c.sh->bar, c.phase, c.err)) c.sh->abort = 1;
  c.phase ^= 1;
  __syncthreads();
  return !c.sh->abort;
}

// x 2^e for |e| <= 126 by one exact multiplication, else ldexpf.
GLA_DEV float scale2(float x, int e) {
  return (e >= -126 && e <= 126) ? x * __int_as_float((e + 127) << 23) : ldexpf(x, e);
}

// Seven slices of the pair (v0, v1) / 2^e into dst + s * stride (bf16x2),
// as k_oz_tile: d = rint(128 v), then the remainder times 128, kept exactly
// in double-float. th - d is a multiple of ulp(th) and |tl| <= ulp(th) / 2,
// so the remainder's (hi, lo) comes from a fast two-sum.
GLA_DEV void slice7x2(df64 v0, df64 v1, int e, unsigned char* dst, int stride) {
  float h0 = scale2(v0.hi, -e), l0 = scale2(v0.lo, -e);
  float h1 = scale2(v1.hi, -e), l1 = scale2(v1.lo, -e);
#pragma unroll
  for (int s = 0; s < kS; s++) {
    const float t0 = h0 * 128.f, u0 = l0 * 128.f, t1 = h1 * 128.f, u1 = l1 * 128.f;
    const float d0 = rintf(t0), d1 = rintf(t1);
    quick_two_sum(t0 - d0, u0, h0, l0);
    quick_two_sum(t1 - d1, u1, h1, l1);
    *reinterpret_cast<__nv_bfloat162*>(dst + s * stride) = __floats2bfloat162_rn(d0, d1);
  }
}

GLA_DEV int exp_of(float m) { return m > 0.f ? ilogbf(m) + 1 : 0; }

// Scale exponents of the columns of an n x n column-major array: out[j] =
// exp_of(max_k |hi(M(k, j))|), one warp per column, four columns in flight
// per warp (all threads of the CTA; ends with a barrier). A row of P whose
// exponent is given this way (P = X', or P = A symmetric) needs no pass of
// its own.
template <class T>
GLA_DEV float hi_of(const T& v);
template <>
GLA_DEV float hi_of<float>(const float& v) { return v; }
template <>
GLA_DEV float hi_of<df64>(const df64& v) { return v.hi; }
template <class T>
GLA_DEV void col_exps(int n, const T* __restrict__ M, int* out) {
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int j0 = wid * 4; j0 < n; j0 += nw * 4) {
    float m[4] = {0.f, 0.f, 0.f, 0.f};
    for (int k = lane; k < n; k += 32)
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (j0 + u < n) m[u] = fmaxf(m[u], fabsf(hi_of(M[(size_t)(j0 + u) * n + k])));
#pragma unroll
    for (int u = 0; u < 4; u++) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) m[u] = fmaxf(m[u], __shfl_xor_sync(0xffffffffu, m[u], o));
      if (lane == 0 && j0 + u < n) out[j0 + u] = exp_of(m[u]);
    }
  }
  __syncthreads();
}

// Scale exponents of the rows of an n x n column-major array: out[i] =
// exp_of(max_j |hi(M(i, j))|), one thread per row (consecutive threads read
// consecutive rows of a column); all threads of the CTA, ends with a barrier.
template <class T>
GLA_DEV void row_exps(int n, const T* __restrict__ M, int* out) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    float m = 0.f;
#pragma unroll 4
    for (int j = 0; j < n; j++) m = fmaxf(m, fabsf(hi_of(M[(size_t)j * n + i])));
    out[i] = exp_of(m);
  }
  __syncthreads();
}

// Slab staging: a warp fills whole 8 x 8 core matrices (each lane one row
// and two consecutive k: 128 contiguous bytes per warp and slice, free of
// bank conflicts). P's 128 x 32 slab is 64 core matrices (8 per warp), Q's
// 32 x 32 slab 16 (2 per warp). The values are loaded into registers first
// (all loads of a slab in flight together) and sliced after.
constexpr int kPPairs = kM * kKS / 2 / 256;   // pairs per thread: 8
constexpr int kQPairs = kNT * kKS / 2 / 256;  // 2
struct SlabRegs {
  df64 p[kPPairs][2];
  df64 q[kQPairs][2];
};

// core matrix cm of a slab with rows/8 row groups: rows 8 (cm / 4) + lane / 4,
// k 8 (cm % 4) + 2 (lane % 4)
GLA_DEV int cm_row(int cm, int lane) { return ((cm >> 2) << 3) + (lane >> 2); }
GLA_DEV int cm_k(int cm, int lane) { return ((cm & 3) << 3) + ((lane & 3) << 1); }

// rows: the rows of P this pass needs (the rest are zero slices); nc: the
// columns of Q.
template <class LP, class LQ>
GLA_DEV void slab_load(SlabRegs& g, int n, int nc, int rows, int k0, int j0, const LP& lp, const LQ& lq) {
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const df64 zero = df_make(0.f, 0.f);
#pragma unroll
  for (int t = 0; t < kPPairs; t++) {
    const int cm = wid + 8 * t;
    const int r = cm_row(cm, lane), k = k0 + cm_k(cm, lane);
    g.p[t][0] = (r < rows && k < n) ? lp(r, k) : zero;
    g.p[t][1] = (r < rows && k + 1 < n) ? lp(r, k + 1) : zero;
  }
#pragma unroll
  for (int t = 0; t < kQPairs; t++) {
    const int cm = wid + 8 * t;
    const int j = j0 + cm_row(cm, lane), k = k0 + cm_k(cm, lane);
    g.q[t][0] = (j < nc && k < n) ? lq(k, j) : zero;
    g.q[t][1] = (j < nc && k + 1 < n) ? lq(k + 1, j) : zero;
  }
}

// doP = false: Q's slab only (P's comes from the cache).
GLA_DEV void slab_slice(const SlabRegs& g, const Ctx& c, int nc, int rows, int j0, const int* ea, const int* eb,
                        bool doP) {
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* sa = c.slabs;
  unsigned char* sb = c.slabs + kS * kABlk;
#pragma unroll
  for (int t = 0; t < kPPairs; t++) {
    if (!doP) break;
    const int cm = wid + 8 * t;
    const int r = cm_row(cm, lane), kk = cm_k(cm, lane);
    unsigned char* dst = sa + oz::tile_off(r, kk);
    if (r < rows) {
      slice7x2(g.p[t][0], g.p[t][1], ea[r], dst, kABlk);
    } else {  // rows of the M = 128 operand not needed (or beyond n)
#pragma unroll
      for (int q = 0; q < kS; q++) *reinterpret_cast<uint32_t*>(dst + q * kABlk) = 0u;
    }
  }
#pragma unroll
  for (int t = 0; t < kQPairs; t++) {
    const int cm = wid + 8 * t;
    const int cc = cm_row(cm, lane), kk = cm_k(cm, lane);
    const int j = j0 + cc;
    unsigned char* dst = sb + oz::tile_off(cc, kk);
    if (j < nc) {
      slice7x2(g.q[t][0], g.q[t][1], eb[j], dst, kBBlk);
    } else {
#pragma unroll
      for (int q = 0; q < kS; q++) *reinterpret_cast<uint32_t*>(dst + q * kBBlk) = 0u;
    }
  }
}

// C = P Q for n <= 128 (all 256 threads of the CTA). ea[i] / eb[j]: scale
// exponents of row i of P and column j of Q (shared memory, i, j < n; any
// e with 2^e >= the row's or column's largest |hi| is exact, the smallest
// such is the most accurate). upper: only i <= j is stored. Returns false
// when the CTA has aborted (C is then incomplete).
template <class LP, class LQ, class ST>
GLA_DEV bool gemm(Ctx& c, int n, int nc, const int* ea, const int* eb, const LP& lp, const LQ& lq, const ST& store,
                  bool upper) {
  const int tid = threadIdx.x;
  if (c.sh->abort) return false;
  const int nks = (n + kKS - 1) / kKS;
  // the P cache pays from the second pass on (n > 32)
  const bool cache = c.pcache != nullptr && nc > kNT;
  SlabRegs g;
  for (int j0 = 0; j0 < nc; j0 += kNT) {
    const bool from_cache = cache && j0 > 0;
    // P rows sliced: all; or (upper, no cache) the stored i <= j < j0 + 32
    const int rows = (upper && !cache) ? min(n, j0 + kNT) : n;
    slab_load(g, n, nc, from_cache ? 0 : rows, 0, j0, lp, lq);
    if (from_cache && j0 == kNT && tid == 0) bulk_wait_all();  // pass 0's stores have landed
    for (int q = 0; q < nks; q++) {
      // the MMAs of the previous slab read the buffers (and, in pass 0 with
      // the cache, its bulk store read P's part): wait for them
      if (q > 0) {
        if (cache && !from_cache && tid == 0) bulk_wait_read();
        if (!wait_mma(c)) return false;
      }
      if (from_cache) {
        if (tid == 0) {
          c.sh->ld_pending = 1;
          c.sh->ld_parity = c.ldphase;
          oz::mbar_expect_tx(&c.sh->ldbar, (uint32_t)kPSlab);
          oz::bulk_g2s(c.slabs, c.pcache + (size_t)q * kPSlab, (uint32_t)kPSlab, &c.sh->ldbar);
        }
        slab_slice(g, c, nc, rows, j0, ea, eb, false);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const bool landed = oz::mbar_wait(&c.sh->ldbar, c.ldphase, c.err);
        c.ldphase ^= 1;
        if (!landed) c.sh->abort = 1;
        __syncthreads();
        if (c.sh->abort) return false;
        if (tid == 0) c.sh->ld_pending = 0;
      } else {
        slab_slice(g, c, nc, rows, j0, ea, eb, true);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
      }
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint64_t a0 = oz::make_desc(oz::smem_u32(c.slabs));
        const uint64_t b0 = oz::make_desc(oz::smem_u32(c.slabs + kS * kABlk));
#pragma unroll
        for (int ks = 0; ks < kKS / 16; ks++)
#pragma unroll
          for (int s = 1; s <= kS; s++) {
            // slice s of P times slices 1 .. 8 - s of Q into levels s + 1 .. 8;
            // s = 1 reaches every level first, so its MMA of the pass's first
            // k step starts the accumulators from zero
            const uint32_t acc = (q == 0 && ks == 0 && s == 1) ? 0u : 1u;
            oz::mma_f16(c.sh->tmem + (uint32_t)((s - 1) * kNT), a0 + (uint64_t)(((s - 1) * kABlk + ks * 256) >> 4),
                        b0 + (uint64_t)((ks * 256) >> 4), idesc_n(kNT * (kS + 1 - s)), acc);
          }
        oz::mma_commit(&c.sh->bar);
        if (cache && !from_cache) bulk_s2g(c.pcache + (size_t)q * kPSlab, c.slabs, (uint32_t)kPSlab);
      }
      // the next slab's loads overlap these MMAs
      if (q + 1 < nks) slab_load(g, n, nc, from_cache ? 0 : rows, (q + 1) * kKS, j0, lp, lq);
    }
    if (!wait_mma(c)) return false;
    asm volatile("tcgen05.fence::after_thread_sync;");
    // drain: TMEM lane = row of C
    {
      const int wid = tid >> 5, lane = tid & 31;
      const int quarter = wid & 3, half = wid >> 2;
      const int r = quarter * 32 + lane;
      float ph[16], pl[16];
#pragma unroll
      for (int u = 0; u < 16; u++) ph[u] = pl[u] = 0.f;
#pragma unroll 1
      for (int L = kS + 1; L >= 2; L--) {
        uint32_t v[16];
        oz::tmem_ld16(c.sh->tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)((L - 2) * kNT + half * 16), v);
        asm volatile("tcgen05.wait::ld.sync.aligned;");
        const float sc = __int_as_float((127 - 7 * L) << 23);  // 2^(-7 L), L <= 8
#pragma unroll
        for (int u = 0; u < 16; u++) {
          float sh, se;
          two_sum(ph[u], __uint_as_float(v[u]) * sc, sh, se);
          ph[u] = sh;
          pl[u] += se;
        }
      }
      if (r < n) {
        const int er = ea[r];
#pragma unroll
        for (int u = 0; u < 16; u++) {
          const int j = j0 + half * 16 + u;
          if (j >= nc || (upper && r > j)) continue;
          float ah, al;
          two_sum(ph[u], pl[u], ah, al);
          const int e = er + eb[j];
          store(r, j, df_make(scale2(ah, e), scale2(al, e)));
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();  // the accumulators are free for the next pass
  }
  return true;
}

// C = P Q with Q square (nc = n).
template <class LP, class LQ, class ST>
GLA_DEV bool gemm(Ctx& c, int n, const int* ea, const int* eb, const LP& lp, const LQ& lq, const ST& store,
                  bool upper) {
  return gemm(c, n, n, ea, eb, lp, lq, store, upper);
}

}  // namespace tcs
}  // namespace gla
