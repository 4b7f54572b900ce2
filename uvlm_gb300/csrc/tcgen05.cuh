// Blackwell (sm_100a / sm_103a) tensor-core primitives in inline PTX:
// tensor memory (TMEM) allocation, tcgen05.mma with the A operand in TMEM and
// the B operand in shared memory, tcgen05.commit to an mbarrier, TMEM
// loads/stores, the tcgen05 ordering fences, and bounded mbarrier waits.
//
// Layouts used here (single CTA, cta_group::1):
//  * D (accumulator, FP32) and A (M x K, one 32-bit element per column):
//    TMEM lane = row, TMEM column = column / K index.  Warp w of a 128-thread
//    block reads and writes lanes 32w .. 32w + 31 (its quarter of TMEM).
//  * B (K x N), K-major without swizzle: built from 8 x 16-byte core
//    matrices (8 consecutive N rows, 16 bytes of K each); the descriptor's
//    leading byte offset is the distance between core matrices adjacent in
//    K, its stride byte offset the distance between core matrices adjacent
//    in N.
#pragma once
#include <cstdint>

namespace vfmm {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ---- tensor memory ----------------------------------------------------------
// Allocate `ncols` TMEM columns (power of two, >= 32); the base address is
// written to shared memory at `dst`.  Executed by one whole warp.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() { asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// TMEM address of lane `lane` and column `col` relative to `base`.
__device__ __forceinline__ uint32_t tmem_addr(uint32_t base, int lane, int col) { return base + ((uint32_t)lane << 16) + (uint32_t)col; }

// 32 lanes x 32 bits, 8 consecutive columns per thread (thread t of the warp:
// lane base + t).
__device__ __forceinline__ void tmem_st8(uint32_t taddr, const uint32_t (&v)[8])
{
  asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr), "r"(v[0]), "r"(v[1]), "r"(v[2]),
               "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7])
               : "memory");
}
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, uint32_t (&v)[8])
{
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7])
               : "r"(taddr)
               : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---- ordering -----------------------------------------------------------------
// tcgen05 operations before a thread barrier / after it.
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Shared-memory writes of this thread (generic proxy) visible to the tensor
// core's reads (async proxy).
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// x rounded to the nearest TF32 value (ties away from zero), as an FP32 bit
// pattern with the 13 low mantissa bits zero; x - tf32_rn(x) is exact in FP32.
__device__ __forceinline__ float tf32_rn(float v)
{
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(v));
  return __uint_as_float(r & 0xFFFFE000u);
}

// ---- descriptors --------------------------------------------------------------
// Shared-memory matrix descriptor, no swizzle: start address, leading byte
// offset (K direction), stride byte offset (M/N direction); bit 46 is the
// fixed descriptor version of sm_100.
__device__ __forceinline__ uint64_t smem_desc_noswizzle(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
         (1ull << 46);
}
// Instruction descriptor of kind::tf32: D FP32, A and B TF32, both K-major,
// no negation, M x N.
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N)
{
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---- MMA ----------------------------------------------------------------------
// D (TMEM) = A (TMEM) x B (shared memory) [+ D if accumulate]; one thread issues.
__device__ __forceinline__ void mma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc, uint32_t accumulate)
{
  asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
               "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
               "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
               : "memory");
}
// Arrive once on `mbar` when every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint64_t *mbar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// ---- mbarrier -----------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *b, uint32_t parity)
{
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok)
               : "r"(smem_u32(b)), "r"(parity)
               : "memory");
  return ok != 0;
}
// Wait for the phase with `parity` to complete, for at most ~`limit` clock
// cycles; false when the limit ran out (the caller records an error).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *b, uint32_t parity, long long limit = 2000000000ll)
{
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity))
    if (clock64() - t0 > limit)
      return false;
  return true;
}

} // namespace tc
} // namespace vfmm
