// tcgen05 building blocks shared by the tensor-core Ozaki GEMMs: the
// canonical no-swizzle K-major shared-memory layout of bf16 operand slabs,
// its matrix descriptor, bounded mbarrier waits, bulk copies, the MMA issue
// and commit, TMEM loads, and the scale exponent of a slice set.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "gla_common.cuh"

namespace gla {
namespace oz {

constexpr int kKS = 32;  // k per slab (two K = 16 MMAs per slice pair)
constexpr long long kWaitLimit = 1ll << 26;

// Byte offset of element (r, kk) inside a tiled slab block (8-row x 8-k core
// matrices of 128 contiguous bytes; K-neighbours 128 B apart = LBO, row
// groups kSBO = 512 B apart = SBO).
constexpr int kSBO = kKS * 16;
__host__ __device__ __forceinline__ int tile_off(int r, int kk) {
  return (r >> 3) * kSBO + (kk >> 3) * 128 + (r & 7) * 16 + (kk & 7) * 2;
}

GLA_DEV uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

GLA_DEV uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;  // LBO: K-neighbour core matrices
  d |= (uint64_t)(((uint32_t)kSBO >> 4) & 0x3FFF) << 32;  // SBO: next 8-row group
  d |= (uint64_t)1 << 46;                        // descriptor version (tcgen05)
  return d;                                      // base offset 0, no swizzle
}


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
GLA_DEV void mma_f16(uint32_t tmem_d, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\ntcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(
          tmem_d),
      "l"(ad), "l"(bd), "r"(idesc), "r"(accumulate));
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

GLA_DEV int slice_exp(unsigned mb) {
  const float m = __uint_as_float(mb);
  return m > 0.f ? ilogbf(m) + 1 : 0;
}

}  // namespace oz
}  // namespace gla
