// grid_sync.cuh — grid-wide barrier of a cooperative launch (device).
#pragma once

#include <cstdint>

#include "world.h"

namespace axiom_gb300 {

constexpr uint32_t kErrBarrier = 8u;  // DevCounters::errorFlags: a grid-barrier wait gave up
constexpr uint32_t kBarrierSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t ldAcquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Every CTA's thread 0 arrives on a monotonic counter and waits for `target` arrivals
// (all CTAs of a cooperative launch are resident, so every wait ends).  The wait is still
// bounded: past the limit, or once another CTA has given up, it sets kErrBarrier and
// returns false, and the caller leaves the kernel instead of hanging.
__device__ __forceinline__ bool gridBarrier(uint32_t* bar, uint32_t target, DevCounters* cnt) {
    __shared__ uint32_t ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(bar, 1u);
        uint32_t it = 0;
        uint32_t good = 1u;
        while (ldAcquire(bar) < target) {
            if (++it > kBarrierSpinLimit || (it % 1024u == 0u && (ldAcquire(&cnt->errorFlags) & kErrBarrier))) {
                atomicOr(&cnt->errorFlags, kErrBarrier);
                good = 0u;
                break;
            }
            __nanosleep(32);
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0u;
}

}  // namespace axiom_gb300
