// tcgen05.cuh — thin inline-PTX wrappers for the 5th-generation tensor core (sm_103a).
//
// Operands live in shared memory in the K-major, no-swizzle canonical layout: "core
// matrices" of 8 rows x 16 bytes (8 bf16 along K) stored contiguously (128 B).  A tile of
// R rows x 64 K-elements puts core matrix (row group g, K chunk c) at byte
// (g * 8 + c) * 128, so the K-direction core-matrix stride (LBO) is 128 B and the 8-row
// group stride (SBO) is 1024 B.  One MMA (kind::f16, K = 16) covers two K chunks; the
// next MMA starts 256 B further.  The fp32 accumulator lives in tensor memory: row i of
// the M = 128 tile is TMEM lane i, column j is TMEM column base + j.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace axiom_gb300 {
namespace tc {

__device__ __forceinline__ uint32_t smemAddr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05): start, leading and stride byte offsets in
// 16-byte units, descriptor version 1, base offset 0, no swizzle.
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;  // version
    return d;                 // layout type 0 (no swizzle) in bits 61-63
}

// Instruction descriptor, kind::f16: BF16 x BF16 -> F32, both operands K-major.
__host__ __device__ constexpr uint32_t idescBf16F32(uint32_t m, uint32_t n) {
    return (1u << 4)            // D format F32
           | (1u << 7)          // A format BF16
           | (1u << 10)         // B format BF16
           | ((n >> 3) << 17)   // N / 8
           | ((m >> 4) << 24);  // M / 16
}

// Warp-wide: allocate ncols TMEM columns, address written to *dst (shared memory).
__device__ __forceinline__ void tmemAlloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smemAddr(dst)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
}

__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
// Makes generic-proxy shared-memory writes visible to the tensor core (async proxy).
__device__ __forceinline__ void fenceProxyAsync() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// Single thread: D (+)= A * B^T, one K = 16 step.
__device__ __forceinline__ void mmaBf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Single thread: arrive on the mbarrier when all prior tcgen05.mma of this thread finish.
__device__ __forceinline__ void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                     smemAddr(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbarInit(uint64_t* mbar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smemAddr(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

// Bounded wait for the phase with the given parity; false after maxSpins polls.
__device__ __forceinline__ bool mbarWait(uint64_t* mbar, uint32_t parity, uint32_t maxSpins) {
    const uint32_t a = smemAddr(mbar);
    for (uint32_t i = 0; i < maxSpins; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Warp-wide: 32 lanes x 16 consecutive fp32 columns of TMEM into v[0..15].
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of element (row, k) of a K-major no-swizzle tile whose K chunk is 64 wide.
__host__ __device__ constexpr uint32_t coreOffset(uint32_t row, uint32_t k) {
    return (((row >> 3) * 8u + (k >> 3)) * 128u) + ((row & 7u) * 16u) + ((k & 7u) * 2u);
}

}  // namespace tc
}  // namespace axiom_gb300
