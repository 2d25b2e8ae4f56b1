// Blackwell (sm_103a) tensor-core primitives for the warm-start network:
// tcgen05 MMA with accumulators in tensor memory (TMEM), operands staged in
// shared memory by TMA tensor copies, completion tracked by mbarriers.
//
// Operand layouts are the tcgen05 "canonical" shared-memory layouts with the
// 64-byte swizzle: rows of 64 bytes (32 bf16), eight-row groups 512 bytes
// apart, 16-byte chunks of row r XOR-permuted by (r >> 1) & 3 -- exactly what
// a TMA tiled copy with CU_TENSOR_MAP_SWIZZLE_64B writes for a box whose
// inner extent is 32 bf16.  Every staged tile starts on a 1024-byte boundary.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace opyx {
namespace tc {

// Iteration bound of every mbarrier wait (each try_wait may itself suspend
// for a while); on expiry the waiting role records a fault and leaves.
constexpr unsigned kSpin = 1u << 22;

OPYX_D uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

OPYX_D void mbar_init(uint64_t* m, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}

OPYX_D void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

OPYX_D void mbar_expect_tx(uint64_t* m, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes)
               : "memory");
}

OPYX_D bool mbar_try(uint64_t* m, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(m)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.
OPYX_D bool mbar_wait(uint64_t* m, unsigned parity) {
  for (unsigned i = 0; i < kSpin; ++i)
    if (mbar_try(m, parity)) return true;
  return false;
}

// TMA tiled loads (global -> shared), completing on an mbarrier.
OPYX_D void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* m) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(m))
      : "memory");
}

OPYX_D void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                        uint64_t* m) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(m))
      : "memory");
}

OPYX_D void prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)map) : "memory");
}

// ---- tensor memory
// Warp-wide: allocates `ncols` (a power of two >= 32) columns x 128 lanes
// and writes the base address to *dst.
OPYX_D void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
               "r"(ncols)
               : "memory");
}
OPYX_D void tmem_relinquish() {
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
OPYX_D void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
OPYX_D void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
OPYX_D void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- descriptors
// Instruction descriptor of kind::f16 with BF16 A and B, FP32 accumulator,
// both operands K-major (a_mn / b_mn select MN-major), M x N tile.
OPYX_HD uint32_t idesc_bf16(int M, int N, int a_mn = 0, int b_mn = 0) {
  return (1u << 4)                      // D format: F32
         | (1u << 7)                    // A format: BF16
         | (1u << 10)                   // B format: BF16
         | ((uint32_t)a_mn << 15)       // A major-ness
         | ((uint32_t)b_mn << 16)       // B major-ness
         | ((uint32_t)(N >> 3) << 17)   // N / 8
         | ((uint32_t)(M >> 4) << 24);  // M / 16
}

// Shared-memory matrix descriptor, 64-byte swizzle.  lbo / sbo in bytes:
// K-major: sbo = stride of eight-row groups (512 for packed 64-byte rows),
// lbo unused; MN-major: lbo = stride between 32-element blocks along M/N,
// sbo = stride of eight-row groups along K.
OPYX_D uint64_t sdesc_sw64(const void* smem, uint32_t lbo, uint32_t sbo) {
  const uint32_t a = smem_u32(smem);
  return (uint64_t)((a >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46)  // descriptor version (sm_100 family)
         | (4ull << 61);                                           // layout: 64-byte swizzle
}

// D[tmem] (+)= A * B^T over one K = 16 slice (kind::f16, one CTA).
OPYX_D void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)acc)
      : "memory");
}

// Arrive on `m` once every MMA issued so far by this thread has completed.
OPYX_D void mma_commit(uint64_t* m) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_u32(m))
               : "memory");
}

// 32 lanes x 16 columns of 32-bit accumulator: thread t of the warp gets
// lane (taddr lane + t), columns [col, col + 16).
OPYX_D void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
}
OPYX_D void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

}  // namespace tc
}  // namespace opyx
