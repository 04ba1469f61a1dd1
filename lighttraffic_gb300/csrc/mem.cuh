// mem.cuh -- loads and reductions with L2 eviction-priority hints.
//
// A random walk reads three streams per hop: the row offsets of the current
// vertex, one column entry, and (PageRank) one counter.  Column entries are
// scattered over the whole col array and are almost never reused, while the
// row offsets and counters of hub vertices are reused constantly.  Marking
// the column loads evict-first (and not allocating them in L1) and the row
// offsets and counters evict-last keeps the reused lines in the 126 MB L2
// instead of letting the column stream flush them.
#pragma once

#include <cstdint>

namespace lt {

__device__ __forceinline__ uint64_t l2_policy_evict_first()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint64_t l2_policy_evict_last()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

// Read-only load through the non-coherent path with an L2 policy.
__device__ __forceinline__ uint64_t ld_nc_u64(const void *a, uint64_t pol)
{
    uint64_t v;
    asm volatile("ld.global.nc.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(a), "l"(pol));
    return v;
}

__device__ __forceinline__ uint32_t ld_nc_u32(const void *a, uint64_t pol)
{
    uint32_t v;
    asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}

// Read-only streaming load: not kept in L1, L2 policy as given.
__device__ __forceinline__ uint32_t ld_nc_stream_u32(const void *a, uint64_t pol)
{
    uint32_t v;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}

// counts[i] += 1 without a return value, with an L2 policy.
__device__ __forceinline__ void red_add1_u64(unsigned long long *a, uint64_t pol)
{
    asm volatile("red.global.add.L2::cache_hint.u64 [%0], 1, %1;" ::"l"(a), "l"(pol) : "memory");
}

// counts[i] += 1 on a u32 counter, with an L2 policy.
__device__ __forceinline__ void red_add1_u32(unsigned int *a, uint64_t pol)
{
    asm volatile("red.global.add.L2::cache_hint.u32 [%0], 1, %1;" ::"l"(a), "l"(pol) : "memory");
}

}  // namespace lt
