// TMA (cp.async.bulk.tensor) and mbarrier helpers for sm_103a, in inline PTX.
//
// Every wait is bounded: bounded_wait() gives up after kWaitLimitNs of
// %globaltimer time and reports false, so a kernel can record an error
// status and return instead of hanging the GPU.  Waiting threads are
// suspended by the hardware (try_wait with a suspend-time hint) instead of
// spinning, so they do not take issue slots from the threads that compute.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace scafes {

// 2 s: far beyond any legitimate TMA latency, short enough to fail fast.
constexpr uint64_t kWaitLimitNs = 2000000000ull;
// Upper bound of one hardware suspension inside try_wait.
constexpr uint32_t kSuspendHintNs = 100000u;

__device__ __forceinline__ uint64_t global_timer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's prior generic-proxy shared-memory accesses before
// subsequent async-proxy (TMA) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// try_wait that lets the hardware suspend the thread for up to `hint_ns`
// while the phase is incomplete.
__device__ __forceinline__ bool mbar_try_wait_suspend(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
        : "memory");
    return ok != 0;
}

// Waits for phase `parity` of `bar` to complete; false once kWaitLimitNs
// (or `limit_ns`) of wall time passed without completion.
__device__ __forceinline__ bool bounded_wait(uint64_t* bar, uint32_t parity,
                                             uint64_t limit_ns = kWaitLimitNs) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_timer_ns();
    while (true) {
        if (mbar_try_wait_suspend(bar, parity, kSuspendHintNs)) return true;
        if (global_timer_ns() - t0 > limit_ns) return false;
    }
}

// 3D tiled TMA load of the box at (x, y, z) into shared memory; completion
// is signalled on `bar` (complete_tx).  x * element size must be a multiple
// of 16 bytes; x, y, z may be negative or beyond the extent (zero fill).
__device__ __forceinline__ void tma_load_3d(void* smem_dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// Host: encodes a 3D tiled tensor map over a padded field
// (dims nx, ny, nz; row pitch and plane pitch in bytes) with box
// (bx, by, 1) elements of `esz` bytes.  Returns CUDA_SUCCESS or the error.
CUresult make_tensor_map_3d(CUtensorMap* map, const void* base, int esz, int nx, int ny, int nz,
                            size_t row_bytes, size_t plane_bytes, int bx, int by);

}  // namespace scafes
