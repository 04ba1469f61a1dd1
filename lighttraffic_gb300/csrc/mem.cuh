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

__device__ __forceinline__ uint2 ld_nc_u2(const void *a, uint64_t pol)
{
    uint2 v;
    asm volatile("ld.global.nc.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(v.x), "=r"(v.y) : "l"(a), "l"(pol));
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

// ---- bulk copies global -> shared (the TMA unit's untiled mode) and the
// mbarriers that count their bytes.  Both addresses and the size must be
// multiples of 16 bytes.

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *m, uint32_t arrivals)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(m)), "r"(arrivals) : "memory");
}

// Makes initialised mbarriers visible to the bulk-copy (async) proxy.
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// One arrival that also announces `bytes` of bulk copies completing on m.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *m, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(m)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *m, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(m)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for the phase of parity `parity` of m to complete; false once
// `limit_ns` have passed (or 2^26 polls) without it.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *m, uint32_t parity, uint64_t limit_ns)
{
    if (mbar_try_wait(m, parity)) return true;
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t k = 0; k < (1u << 26); k++) {
        if (mbar_try_wait(m, parity)) return true;
        if ((k & 63) == 63 && globaltimer_ns() - t0 > limit_ns) return false;
    }
    return false;
}

// Bulk copy of `bytes` from global memory into this CTA's shared memory;
// completion is counted on m.
__device__ __forceinline__ void bulk_load_smem(void *dst, const void *src, uint32_t bytes, uint64_t *m)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"((uint64_t)__cvta_generic_to_global(src)), "r"(bytes), "r"(smem_addr(m))
                 : "memory");
}

}  // namespace lt
