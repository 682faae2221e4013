// tma.cuh -- Tensor Memory Accelerator loads and mbarrier waits (sm_90+ PTX,
// used on sm_103a).  Every wait is bounded: after kTmaSpinLimit polls the
// caller gets false and must set an error flag and leave.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace fp {

constexpr long long kTmaSpinLimit = 1LL << 22;  // polls (each try_wait may sleep briefly)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make the barrier initialisation visible to the async (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// order earlier generic-proxy shared-memory accesses before later async-proxy ones
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase with the given parity to complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (long long it = 0; it < kTmaSpinLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// Acquire fence for a tensor map that lives in global memory (copied there by
// the host before the launch): later TMA copies through it see its contents,
// not a stale copy of an earlier map at the same address.
__device__ __forceinline__ void fence_tensormap_acquire(const CUtensorMap* map) {
    asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(
                     reinterpret_cast<uint64_t>(map))
                 : "memory");
}

// 4-D tiled TMA load global -> shared, completing on bar (transaction bytes).
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
                                            int c3, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// 1-D bulk copy global -> shared, completing on bar (transaction bytes).
// dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// Wait of a two-stage pipeline for stage b of iteration i (parity (i >> 1) & 1).
// Every thread of the CTA calls it.  On a timeout the CTA raises *err, thread 0
// waits (bounded) for its own prefetch of the other stage when one was issued,
// and all threads get false and must return.
template <typename T2>
__device__ __forceinline__ bool tma_pipeline_wait(uint64_t* bars, int i, int b, bool prefetched,
                                                  int* err) {
    const bool ok = mbar_wait_bounded(&bars[b], (uint32_t)((i >> 1) & 1));
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            if (prefetched) mbar_wait_bounded(&bars[b ^ 1], (uint32_t)(((i + 1) >> 1) & 1));
        }
        return false;
    }
    return true;
}

}  // namespace fp
