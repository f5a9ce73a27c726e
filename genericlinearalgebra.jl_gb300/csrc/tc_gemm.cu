// 3xTF32 tcgen05 GEMM with TMA-fed operands (declarations and the numerics
// in tc_gemm.cuh).
//
// CTA: one 128 x 128 tile of D, 256 threads, a 3-stage ring of 64 KB
// stages (A and B tiles of 128 rows x 32 k as loaded, plus their low parts).
//   warp 0 (one lane): TMA loads of A and B into a stage
//     (cp.async.bulk.tensor.2d, 128-byte swizzle, completion on the stage's
//     "full" mbarrier);
//   warps 4-7 (128 threads): split the stage in place, hi = x rounded to TF32,
//     lo = x - hi rounded to TF32 into the stage's low-part tiles (same
//     swizzled offsets), then a proxy fence and an arrive on "split";
//   warp 1 (one lane): per stage 4 k-steps x 3 tcgen05.mma kind::tf32
//     (hi hi, hi lo, lo hi; M = N = 128, K = 8) into one TMEM accumulator of
//     128 columns, then tcgen05.commit to the stage's "empty" mbarrier;
//   all eight warps: after the last commit, tcgen05.ld of the accumulator
//     (each warp a 32-lane quarter = 32 rows of D, and half of the columns)
//     and the alpha/beta store, rows of a column contiguous across the
//     lanes; the first 32 C values of each thread are loaded before the
//     accumulator completes.
// Every mbarrier wait is bounded: a wait that runs out sets the error word
// and the CTA stops issuing work, waits (bounded) for its own copies and
// MMAs, frees its TMEM and returns.
#include <cudaTypedefs.h>

#include <mutex>

#include "../../include/glagpu.h"
#include "gla_common.cuh"
#include "tc_gemm.cuh"

namespace gla {
namespace tc {

namespace {

constexpr int kStages = 3;
constexpr int kTile = kBM * kBK * 4;          // 16 KB (A and B tiles alike: kBN == kBM)
constexpr int kStage = 4 * kTile;             // A hi, B hi, A lo, B lo
constexpr int kSmem = kStages * kStage + 1024;  // + alignment slack
constexpr int kThreads = 256;
constexpr long long kWaitLimit = 1ll << 26;
// kind::tf32 instruction descriptor: F32 accumulate (bits 4-5 = 1), TF32 A
// and B (bits 7-9, 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                            ((uint32_t)(kBM >> 4) << 24);
static_assert(kBN == kBM, "A and B tiles share one size");

GLA_DEV uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory descriptor of a K-major tile in the 128-byte-swizzled
// layout the TMA writes: rows of 128 bytes, 8-row groups 1024 bytes apart
// (SBO), version 1, layout type 2 (128-byte swizzle). The tile starts on a
// 1024-byte boundary; a K offset inside the row adds offset >> 4 to the
// address field.
GLA_DEV uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)(1024 >> 4) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}

GLA_DEV void mbar_init(uint64_t* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count));
}
GLA_DEV bool mbar_try(uint64_t* b, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return done != 0;
}
// Bounded wait; false when it ran out (error word set) or the CTA aborted.
GLA_DEV bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag, int* err) {
  for (long long it = 0; it < kWaitLimit; it++) {
    if (mbar_try(b, parity)) return true;
    if ((it & 1023) == 1023 && *abort_flag) return false;
  }
  atomicExch(err, 1);
  *abort_flag = 1;
  return false;
}
GLA_DEV void mbar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
GLA_DEV void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
GLA_DEV void tma_load(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          su32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(su32(bar))
      : "memory");
}
GLA_DEV void mma_tf32(uint32_t tmem_d, uint64_t ad, uint64_t bd, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(
          tmem_d),
      "l"(ad), "l"(bd), "r"(kIdesc), "r"(accumulate));
}
GLA_DEV void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}
GLA_DEV void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}

// x rounded to the nearest TF32 value (19 bits; ties away from zero):
// exactly representable, so the tensor core reads it unchanged.
GLA_DEV float tf32_rn(float x) { return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u); }

// Split one stage tile in place: hi = tf32(x), lo = tf32(x - hi) (x - hi is
// exact in FP32); x - hi - lo is below 2^-22 |x|.
GLA_DEV void split_tile(float4* hi, float4* lo, int t) {
#pragma unroll 4
  for (int v = t; v < kTile / 16; v += 128) {
    const float4 x = hi[v];
    const float4 h = make_float4(tf32_rn(x.x), tf32_rn(x.y), tf32_rn(x.z), tf32_rn(x.w));
    hi[v] = h;
    lo[v] = make_float4(tf32_rn(x.x - h.x), tf32_rn(x.y - h.y), tf32_rn(x.z - h.z), tf32_rn(x.w - h.w));
  }
}

__global__ void __launch_bounds__(kThreads, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap mA, const __grid_constant__ CUtensorMap mB, const TcArgs g) {
  extern __shared__ unsigned char sm_raw[];
  __shared__ __align__(8) uint64_t full_bar[kStages], split_bar[kStages], empty_bar[kStages], done_bar, fin_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int s_abort_raw;
  volatile int* s_abort = &s_abort_raw;
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(sm_raw) + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int tiles_m = (g.M + kBM - 1) / kBM;
  const int tm = blockIdx.x % tiles_m, tn = blockIdx.x / tiles_m;
  const int row0 = tm * kBM, col0 = tn * kBN;
  if (g.lower && row0 + kBM <= col0) return;  // (uniform) nothing allocated yet
  // K iterations: per segment, or the split's share of the one segment
  int kbeg = 0, kend = g.K[0];
  if (g.ksplit > 0) {
    kbeg = blockIdx.y * g.ksplit;
    kend = min(g.K[0], kbeg + g.ksplit);
  }
  const int it0 = g.ksplit > 0 ? (max(kend - kbeg, 0) + kBK - 1) / kBK : (g.K[0] + kBK - 1) / kBK;
  const int it1 = (g.nseg > 1 && g.ksplit <= 0) ? (g.K[1] + kBK - 1) / kBK : 0;
  const int niter = it0 + it1;
  float* D = g.D + (g.ksplit > 0 ? (long long)blockIdx.y * g.split_stride : 0ll);
  if (tid == 0) {
    for (int i = 0; i < kStages; i++) {
      mbar_init(&full_bar[i], 1);
      mbar_init(&split_bar[i], 128);
      mbar_init(&empty_bar[i], 1);
    }
    mbar_init(&done_bar, 1);
    mbar_init(&fin_bar, 1);
    *s_abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (wid == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_base)),
                 "r"(kBN));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  int* err = g.err;

  if (wid == 0) {
    // ---- producer
    if (lane == 0 && niter > 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mA)) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&mB)) : "memory");
      int issued = 0;
      for (int it = 0; it < niter && !*s_abort; it++) {
        const int st = it % kStages;
        if (it >= kStages && !mbar_wait(&empty_bar[st], ((it / kStages) - 1) & 1, s_abort, err)) break;
        int ax, bx;
        if (it < it0) {
          const int k = (g.ksplit > 0 ? kbeg : 0) + it * kBK;
          ax = g.a_x[0] + k;
          bx = g.b_x[0] + k;
        } else {
          const int k = (it - it0) * kBK;
          ax = g.a_x[1] + k;
          bx = g.b_x[1] + k;
        }
        unsigned char* stg = sm + st * kStage;
        mbar_expect_tx(&full_bar[st], 2 * kTile);
        tma_load(stg, &mA, ax, g.a_y + row0, &full_bar[st]);
        tma_load(stg + kTile, &mB, bx, g.b_y + col0, &full_bar[st]);
        issued = it + 1;
      }
      // the CTA may exit only once its last copies have landed (bounded)
      for (int it = (issued > kStages ? issued - kStages : 0); it < issued; it++)
        for (long long w = 0; w < kWaitLimit && !mbar_try(&full_bar[it % kStages], (it / kStages) & 1); w++) {
        }
    }
  } else if (wid == 1) {
    // ---- MMA issuer
    if (lane == 0 && niter > 0) {
      for (int it = 0; it < niter && !*s_abort; it++) {
        const int st = it % kStages;
        if (!mbar_wait(&split_bar[st], (it / kStages) & 1, s_abort, err)) break;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t base = su32(sm + st * kStage);
        const uint64_t ahi = desc_sw128(base), bhi = desc_sw128(base + kTile);
        const uint64_t alo = desc_sw128(base + 2 * kTile), blo = desc_sw128(base + 3 * kTile);
#pragma unroll
        for (int kk = 0; kk < kBK / 8; kk++) {  // K = 8 per instruction: 32 bytes of each row
          const uint64_t o = (uint64_t)(kk * 32 >> 4);
          mma_tf32(tmem, ahi + o, bhi + o, (it > 0 || kk > 0) ? 1u : 0u);
          mma_tf32(tmem, ahi + o, blo + o, 1u);
          mma_tf32(tmem, alo + o, bhi + o, 1u);
        }
        mma_commit(&empty_bar[st]);
        if (it == niter - 1) mma_commit(&done_bar);
      }
    }
  } else if (wid >= 4) {
    // ---- splitters
    const int t = tid - 128;
    for (int it = 0; it < niter; it++) {
      const int st = it % kStages;
      if (!mbar_wait(&full_bar[st], (it / kStages) & 1, s_abort, err)) break;
      float4* stg = reinterpret_cast<float4*>(sm + st * kStage);
      split_tile(stg, stg + 2 * (kTile / 16), t);                  // A
      split_tile(stg + kTile / 16, stg + 3 * (kTile / 16), t);     // B
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // visible to the tensor core
      mbar_arrive(&split_bar[st]);
    }
  }
  // ---- epilogue, all eight warps: warp w reads TMEM lane quarter w % 4 (rows
  // 32 (w % 4) .. of the tile) and the column half w / 4; the first 32
  // values of C it updates are loaded before the accumulator is complete
  __syncwarp();  // warps 0 and 1 reconverge after their single-lane roles (tcgen05.ld is warp-aligned)
  {
    const int quarter = wid & 3, ch = (wid >> 2) * (kBN / 2);
    const int r = row0 + quarter * 32 + lane;
    const bool rin = r < g.M;
    float cv[32];
    auto load_c = [&](int c0) {
#pragma unroll
      for (int q = 0; q < 32; q++) {
        const int c = col0 + c0 + q;
        cv[q] = 0.f;
        if (g.beta != 0.f && rin && c < g.N && !(g.lower && r < c)) cv[q] = D[(long long)r + (long long)c * g.ldd];
      }
    };
    load_c(ch);
    bool ok = !*s_abort;
    if (ok && niter > 0) ok = mbar_wait(&done_bar, 0, s_abort, err);
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll 1
      for (int c0 = ch; c0 < ch + kBN / 2; c0 += 32) {
        if (c0 != ch) load_c(c0);
        uint32_t v[32];
        if (niter > 0) {
          uint32_t (&v0)[16] = *reinterpret_cast<uint32_t(*)[16]>(&v[0]);
          uint32_t (&v1)[16] = *reinterpret_cast<uint32_t(*)[16]>(&v[16]);
          tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0, v0);
          tmem_ld16(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(c0 + 16), v1);
          asm volatile("tcgen05.wait::ld.sync.aligned;");
        } else {
#pragma unroll
          for (int q = 0; q < 32; q++) v[q] = 0u;
        }
        if (!rin) continue;
#pragma unroll
        for (int q = 0; q < 32; q++) {
          const int c = col0 + c0 + q;
          if (c >= g.N || (g.lower && r < c)) continue;
          D[(long long)r + (long long)c * g.ldd] = fmaf(g.beta, cv[q], g.alpha * __uint_as_float(v[q]));
        }
      }
    }
  }
  // teardown: every MMA of this CTA has finished (a final commit, waited for
  // with a bound) before TMEM is freed
  __syncthreads();
  if (wid == 1 && lane == 0) {
    mma_commit(&fin_bar);
    for (long long w = 0; w < kWaitLimit && !mbar_try(&fin_bar, 0); w++) {
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (wid == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kBN));
}

std::once_flag g_once;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
cudaError_t g_attr = cudaErrorUnknown;

void init_once() {
  std::call_once(g_once, [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &fn, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    g_attr = cudaFuncSetAttribute(k_tc_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
  });
}

}  // namespace

bool tc_available() {
  init_once();
  return g_encode != nullptr && g_attr == cudaSuccess;
}

bool tc_make_map(CUtensorMap* m, const float* base, long long kext, long long rows, long long ld, int box_rows) {
  if (!tc_available()) return false;
  if ((reinterpret_cast<uintptr_t>(base) & 15) != 0 || (ld & 3) != 0 || kext < 1 || rows < 1 || ld < kext)
    return false;
  const cuuint64_t dims[2] = {(cuuint64_t)kext, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box,
                              estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

cudaError_t tc_gemm_launch(const CUtensorMap& mA, const CUtensorMap& mB, const TcArgs& g, int splits,
                           cudaStream_t st) {
  if (g.M <= 0 || g.N <= 0) return cudaSuccess;
  if (!tc_available()) return cudaErrorNotSupported;
  const int tiles = ((g.M + kBM - 1) / kBM) * ((g.N + kBN - 1) / kBN);
  k_tc_gemm<<<dim3(tiles, g.ksplit > 0 ? splits : 1), kThreads, kSmem, st>>>(mA, mB, g);
  return cudaGetLastError();
}

}  // namespace tc
}  // namespace gla

// ---------------------------------------------------------------- C ABI

namespace {
__device__ int g_sgemm_err;  // timeout word of gla_sgemm_3xtf32
std::mutex g_sgemm_mu;
int* g_sgemm_err_addr = nullptr;
}  // namespace

extern "C" int gla_sgemm_3xtf32(int64_t m, int64_t n, int64_t k, float alpha, const float* At, int64_t ldat,
                                const float* B, int64_t ldb, float beta, float* C, int64_t ldc, void* stream) {
  using namespace gla::tc;
  if (m < 0 || m > (1ll << 30)) return -1;
  if (n < 0 || n > (1ll << 30)) return -2;
  if (k < 0 || k > (1ll << 30)) return -3;
  if (!(alpha == alpha)) return -4;
  if ((!At && m && k) || ((uintptr_t)At & 15) != 0) return -5;
  if (ldat < (k > 1 ? k : 1) || (ldat & 3) != 0) return -6;
  if ((!B && n && k) || ((uintptr_t)B & 15) != 0) return -7;
  if (ldb < (k > 1 ? k : 1) || (ldb & 3) != 0) return -8;
  if (!(beta == beta)) return -9;
  if (!C && m && n) return -10;
  if (ldc < (m > 1 ? m : 1)) return -11;
  if (m == 0 || n == 0) return 0;
  if (!tc_available()) return GLA_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_sgemm_mu);
  if (!g_sgemm_err_addr) {
    void* a = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&a, g_sgemm_err);
    if (e != cudaSuccess) return -1000 - (int)e;
    g_sgemm_err_addr = static_cast<int*>(a);
    if ((e = cudaMemset(g_sgemm_err_addr, 0, sizeof(int))) != cudaSuccess) return -1000 - (int)e;
  }
  int h = 0;  // a wait that ran out in an earlier call is reported now
  cudaError_t e = cudaMemcpy(&h, g_sgemm_err_addr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return -1000 - (int)e;
  if (h) {
    cudaMemset(g_sgemm_err_addr, 0, sizeof(int));
    return -1000 - (int)cudaErrorLaunchTimeout;
  }
  CUtensorMap mA, mB;
  if (!tc_make_map(&mA, At, k > 0 ? k : 1, m, ldat, kBM) || !tc_make_map(&mB, B, k > 0 ? k : 1, n, ldb, kBN))
    return GLA_ERR_UNSUPPORTED;
  TcArgs g{};
  g.M = (int)m;
  g.N = (int)n;
  g.nseg = 1;
  g.K[0] = (int)k;
  g.D = C;
  g.ldd = ldc;
  g.alpha = alpha;
  g.beta = beta;
  g.err = g_sgemm_err_addr;
  e = tc_gemm_launch(mA, mB, g, 1, (cudaStream_t)stream);
  return e == cudaSuccess ? 0 : -1000 - (int)e;
}

