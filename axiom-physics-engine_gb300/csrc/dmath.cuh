// dmath.cuh — device fp32 helpers of the rigid-body step.
//
// The whole library is compiled with --fmad=false: every a*b+c below is a rounded
// multiply followed by a rounded add, in the written order, and division and sqrtf are
// IEEE round-to-nearest (nvcc's default -prec-div / -prec-sqrt).  Written that way the
// kernels give bit-identical results to a scalar CPU evaluation of the same expressions.
//
// Semantics follow the reference math layer: Vec3 dot/cross/normalized
// (include/axiom/math/vec3.hpp:179-215), inclusive AABB::intersects
// (include/axiom/math/aabb.hpp:132-135) and the quaternion rotate/normalize of
// src/math/quat.cpp:33-65.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace axd {

struct f3 {
    float x, y, z;
};

__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 mk(float4 v) { return f3{v.x, v.y, v.z}; }
__device__ __forceinline__ f3 add(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 sub(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 scale(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float maxf(float a, float b) { return a > b ? a : b; }
__device__ __forceinline__ float minf(float a, float b) { return a < b ? a : b; }

// v' = (v + w t) + q.xyz x t, t = 2 (q.xyz x v)
__device__ __forceinline__ f3 rotate(float4 q, f3 v) {
    f3 t{2.0f * (q.y * v.z - q.z * v.y), 2.0f * (q.z * v.x - q.x * v.z),
         2.0f * (q.x * v.y - q.y * v.x)};
    return f3{(v.x + q.w * t.x) + (q.y * t.z - q.z * t.y),
              (v.y + q.w * t.y) + (q.z * t.x - q.x * t.z),
              (v.z + q.w * t.z) + (q.x * t.y - q.y * t.x)};
}
__device__ __forceinline__ float4 conj(float4 q) { return make_float4(-q.x, -q.y, -q.z, q.w); }

struct m3 {
    float m[3][3];
};
__device__ __forceinline__ m3 rotmat(float4 q) {
    float xx = q.x * q.x, yy = q.y * q.y, zz = q.z * q.z;
    float xy = q.x * q.y, xz = q.x * q.z, yz = q.y * q.z;
    float wx = q.w * q.x, wy = q.w * q.y, wz = q.w * q.z;
    m3 r;
    r.m[0][0] = 1.0f - 2.0f * (yy + zz);
    r.m[0][1] = 2.0f * (xy - wz);
    r.m[0][2] = 2.0f * (xz + wy);
    r.m[1][0] = 2.0f * (xy + wz);
    r.m[1][1] = 1.0f - 2.0f * (xx + zz);
    r.m[1][2] = 2.0f * (yz - wx);
    r.m[2][0] = 2.0f * (xz - wy);
    r.m[2][1] = 2.0f * (yz + wx);
    r.m[2][2] = 1.0f - 2.0f * (xx + yy);
    return r;
}

// Six unique entries of R diag(i) R^T: (xx, yy, zz, xy), (xz, yz, -, -).
__device__ __forceinline__ float inertiaEntry(const m3& r, f3 i, int a, int b) {
    return r.m[a][0] * i.x * r.m[b][0] + r.m[a][1] * i.y * r.m[b][1] + r.m[a][2] * i.z * r.m[b][2];
}
__device__ __forceinline__ f3 mulSym(float4 s0, float4 s1, f3 v) {
    // s0 = (xx, yy, zz, xy), s1 = (xz, yz, _, _)
    return f3{s0.x * v.x + s0.w * v.y + s1.x * v.z, s0.w * v.x + s0.y * v.y + s1.y * v.z,
              s1.x * v.x + s1.y * v.y + s0.z * v.z};
}

// Duff et al. 2017 orthonormal basis; +0 counts as positive.
__device__ __forceinline__ void tangentBasis(f3 n, f3* t1, f3* t2) {
    float sign = (n.z >= 0.0f) ? 1.0f : -1.0f;
    float a = -1.0f / (sign + n.z);
    float b = n.x * n.y * a;
    *t1 = f3{1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x};
    *t2 = f3{b, sign + n.y * n.y * a, -n.y};
}

__device__ __forceinline__ float4 qnormalize(float4 q) {
    float len = sqrtf(q.x * q.x + q.y * q.y + q.z * q.z + q.w * q.w);
    if (len > 0.0f) {
        float inv = 1.0f / len;
        return make_float4(q.x * inv, q.y * inv, q.z * inv, q.w * inv);
    }
    return q;
}

// SplitMix64 finaliser (a bijection of uint64): colouring priority of a pair key.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t pairKey(uint32_t a, uint32_t b) {
    uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
    return (uint64_t(lo) << 32) | uint64_t(hi);
}

// Block-wide reservation on a global counter: thread i asks for n_i slots and gets the
// first of them; one atomic per block (a counter hit by every warp of a large grid
// serialises in L2).  Every thread of the block calls it; blockDim is a multiple of 32.
__device__ __forceinline__ uint32_t blockReserve(uint32_t n, uint32_t* counter) {
    __shared__ uint32_t warpSum[32];
    __shared__ uint32_t base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = n;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warpSum[warp] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) {
            const uint32_t c = warpSum[w];
            warpSum[w] = total;
            total += c;
        }
        base = total ? atomicAdd(counter, total) : 0u;
    }
    __syncthreads();
    const uint32_t r = base + warpSum[warp] + x - n;
    __syncthreads();  // warpSum / base are reused by the next call
    return r;
}

// Three block-wide reservations in one pass: thread i asks for n0_i, n1_i, n2_i slots (each
// at most 1023 per block in total) on three counters and gets the first of each.  Every
// thread of the block calls it; blockDim is a multiple of 32.
__device__ __forceinline__ uint3 blockReserve3(uint32_t n0, uint32_t n1, uint32_t n2, uint32_t* c0, uint32_t* c1,
                                               uint32_t* c2) {
    __shared__ uint32_t warpSum[32];
    __shared__ uint3 base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t n = n0 | (n1 << 10) | (n2 << 20);
    uint32_t x = n;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) warpSum[warp] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (uint32_t w = 0; w < (blockDim.x >> 5); ++w) {
            const uint32_t c = warpSum[w];
            warpSum[w] = total;
            total += c;
        }
        const uint32_t t0 = total & 1023u, t1 = (total >> 10) & 1023u, t2 = total >> 20;
        base = make_uint3(t0 ? atomicAdd(c0, t0) : 0u, t1 ? atomicAdd(c1, t1) : 0u, t2 ? atomicAdd(c2, t2) : 0u);
    }
    __syncthreads();
    const uint32_t r = warpSum[warp] + x - n;  // this thread's exclusive offsets, packed
    const uint3 b = base;
    __syncthreads();  // warpSum / base are reused by the next call
    return make_uint3(b.x + (r & 1023u), b.y + ((r >> 10) & 1023u), b.z + (r >> 20));
}

}  // namespace axd
