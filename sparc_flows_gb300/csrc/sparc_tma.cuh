// sparc_tma.cuh -- Tensor Memory Accelerator (TMA) and mbarrier helpers (inline PTX, sm_90+).
//
// Tiles of x-fastest fields are moved global -> shared with 2-D tiled bulk tensor copies
// (cp.async.bulk.tensor.2d) completing on a shared-memory mbarrier.  Every wait is bounded: on
// time-out the caller records an error and keeps waiting (again bounded) for the copies it
// issued before leaving, so no copy lands in shared memory of a finished block.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

namespace sparc {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make the initialised barrier visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on phase `parity`; returns false if max_iter polls did not see it complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, uint32_t max_iter)
{
    for (uint32_t i = 0; i < max_iter; i++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 2-D tiled load of box {box_x, box_y} at element coordinates (x, y) into shared memory.
__device__ __forceinline__ void tma_load_2d(void *smem_dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Make this thread's generic-proxy shared-memory accesses visible to / ordered before later
// async-proxy (TMA) operations on the same shared memory.
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// The tensor maps one column pass reads (2-D views [rows][nx] of x-fastest fields).
struct ColMaps {
    CUtensorMap A;    // rows (b*4 + f)*nz + k
    CUtensorMap SV;   // rows ((slot*nb + b)*2 + c)*nz + k
    CUtensorMap DX;   // rows b*nz + k
    CUtensorMap FXX;
    CUtensorMap FXZ;
    CUtensorMap C2R;  // rows b*nz + k (per-solve background) or k (shared)
    CUtensorMap V0Z;  // as C2R
};

// Tensor maps of the 32-column banded column pass (box: 32 columns x nz/2 rows): the state A,
// the RHS ring SV and the row pass's dxi_x/dx, rows as in ColMaps.
struct ColMaps32 {
    CUtensorMap A;
    CUtensorMap SV;
    CUtensorMap DX;  // rows b*nz + k
};

}  // namespace sparc
