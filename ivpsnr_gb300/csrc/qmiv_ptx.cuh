// Inline-PTX helpers for the bulk-copy (TMA) staging: mbarriers and 2-D tensor loads.
#pragma once
#include <cstdint>

namespace qmiv {
namespace ptx {

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\t"
               "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
               "selp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// Bounded wait: gives up after `limit` polls and returns false (the caller records an error).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit)
{
  for(uint32_t i = 0; i < limit; i++)
    if(mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void prefetch_tmap(const void* tmap)
{
  asm volatile("prefetch.tensormap [%0];" :: "l"(tmap) : "memory");
}

// 2-D tiled tensor load into shared memory, completion signalled on `bar` (bytes).
// x must be a multiple of 16 bytes / element size; negative or out-of-range boxes read zeros.
__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, int x, int y, uint64_t* bar)
{
  asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
               :: "r"(smem_addr(dst)), "l"(tmap), "r"(x), "r"(y), "r"(smem_addr(bar)) : "memory");
}

// a*b+c as an integer multiply-add (issued to the FMA pipe rather than the ALU pipe)
__device__ __forceinline__ unsigned mad_u32(unsigned a, unsigned b, unsigned c)
{
  unsigned d;
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(c));
  return d;
}

}  // namespace ptx
}  // namespace qmiv
