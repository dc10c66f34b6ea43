// l2hint.cuh -- global loads and stores of blind-rotation accumulators with an
// L2 evict-last cache policy.
//
// The step-outer schedules write every accumulator back after a step and read
// it again one step later, while each step's bootstrapping-key tile streams
// through L2 once. Under the default policy the key lines push accumulators
// out (the 64-bit kernel wrote its 64 MB of accumulators back to DRAM at every
// step). Accumulator accesses carry a fractional evict_last policy
// (createpolicy + .L2::cache_hint), so L2 evicts the streaming key lines
// before them; key loads keep the default policy. The hint changes where
// lines live in L2, not the values: results are unchanged.
//
// The accesses are volatile asm so that they keep their program order with
// the named barriers and fences around them; loads have no memory clobber, so
// other loads can still be scheduled around them.
#pragma once
#include <cstdint>

namespace fheacc {
namespace dev {

__device__ __forceinline__ uint64_t l2_keep_policy()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint4 ld_keep(const uint4 *a, uint64_t pol)
{
    uint4 v;
    asm volatile("ld.global.cg.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(__cvta_generic_to_global(a)), "l"(pol));
    return v;
}

__device__ __forceinline__ void st_keep(uint4 *a, uint4 v, uint64_t pol)
{
    asm volatile("st.global.cg.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(__cvta_generic_to_global(a)),
                 "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "l"(pol)
                 : "memory");
}

__device__ __forceinline__ uint64_t ld_keep64(const uint64_t *a, uint64_t pol)
{
    uint64_t v;
    asm volatile("ld.global.cg.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(v) : "l"(__cvta_generic_to_global(a)), "l"(pol));
    return v;
}

__device__ __forceinline__ void st_keep64(uint64_t *a, uint64_t v, uint64_t pol)
{
    asm volatile("st.global.cg.L2::cache_hint.u64 [%0], %1, %2;" ::"l"(__cvta_generic_to_global(a)), "l"(v), "l"(pol)
                 : "memory");
}

}  // namespace dev
}  // namespace fheacc
