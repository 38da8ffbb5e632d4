// Shared definitions for the netsci_gb300 CUDA library: status codes, error
// capture, and the small device helpers the KSG and Hedetniemi kernels share.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "errors.h"

// ---------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------

// Chebyshev helpers. Distances are |x_i - x_j| rounded once (subtract) and
// then combined with exact max operations, the arithmetic of
// netcalc/src/mutual_information_cpu.cpp:28-46, so every distance and every
// comparison is bit-identical to the reference CPU path.
__device__ __forceinline__ float nsg_absdiff(float a, float b) { return fabsf(a - b); }

// Three-input maximum (sm_100+ PTX form, one instruction).
__device__ __forceinline__ float nsg_max3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

__device__ __forceinline__ float nsg_min3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Packed pair subtraction: two IEEE round-to-nearest subtractions in one
// instruction on sm_100+ (sub.rn.f32x2); bit-identical to two scalar FSUBs.
// The operands are assembled and split with register-pair moves so no
// extra arithmetic is generated around the packed instruction.
__device__ __forceinline__ void nsg_sub2(float a0, float a1, float b0, float b1, float& r0,
                                         float& r1) {
    asm("{\n\t.reg .b64 pa, pb, pr;\n\t"
        "mov.b64 pa, {%2, %3};\n\t"
        "mov.b64 pb, {%4, %5};\n\t"
        "sub.rn.f32x2 pr, pa, pb;\n\t"
        "mov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r0), "=f"(r1)
        : "f"(a0), "f"(a1), "f"(b0), "f"(b1));
}

__device__ __forceinline__ float2 nsg_sub2(float2 a, float2 b) {
    float2 r;
    nsg_sub2(a.x, a.y, b.x, b.y, r.x, r.y);
    return r;
}

// 1.0f when a <= b, else 0.0f (also when either is NaN): one set.le.f32.f32.
// Counting with these and float adds keeps the count loops off the integer
// select-and-add path (exact while a count stays below 2^24).
__device__ __forceinline__ float nsg_le_f32(float a, float b) {
    float r;
    asm("set.le.f32.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}

// Packed add of two float pairs (add.rn.f32x2), assembled the same way.
__device__ __forceinline__ float2 nsg_add2(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 pa, pb, pr;\n\t"
        "mov.b64 pa, {%2, %3};\n\t"
        "mov.b64 pb, {%4, %5};\n\t"
        "add.rn.f32x2 pr, pa, pb;\n\t"
        "mov.b64 {%0, %1}, pr;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

// Bounded mbarrier wait (phase parity). Returns false when the iteration
// limit runs out; callers record FAULT_WAIT_TIMEOUT and leave.
__device__ __forceinline__ bool nsg_mbar_wait(uint32_t bar_smem, uint32_t parity,
                                              uint32_t max_iters) {
    for (uint32_t it = 0; it < max_iters; ++it) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(bar_smem), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

__device__ __forceinline__ uint32_t nsg_smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// mbarrier and bulk-copy (TMA) primitives.
__device__ __forceinline__ void nsg_mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
// Makes initialised barriers visible to the asynchronous (copy) proxy.
__device__ __forceinline__ void nsg_fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Orders this thread's earlier shared-memory accesses before later
// asynchronous-proxy accesses (a bulk copy into a buffer just read).
__device__ __forceinline__ void nsg_fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
// Arrive on the barrier, announcing `bytes` of asynchronous transfers.
__device__ __forceinline__ void nsg_mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
}
// One-dimensional bulk copy global -> shared, completing on `bar`.
// dst and src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void nsg_bulk_load(uint32_t dst, const void* src, uint32_t bytes,
                                              uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(dst), "l"(src), "r"(bytes), "r"(bar)
        : "memory");
}
